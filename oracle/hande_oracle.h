/*
 * hande_oracle.h -- CPU restatement of HANDE's FCIQMC cycle.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle the GPU engine is checked
 * against: only tests/, __graft_entry__.smoke() and bench.py's CPU baseline
 * load it.  The product library (libhande_gpu.so) never links or calls it.
 *
 * The reference (HANDE, Fortran) cannot be compiled in this environment, so
 * the oracle restates its algorithm function by function, each citing the
 * reference file:line it follows.  It is pinned against the FCI energies of
 * the reference's own test suite (tests/golden/), which fix the Hamiltonian
 * (Slater-Condon rules, integral indexing, k-space symmetry tables).
 *
 * The random numbers come from the same counter-based Philox4x32-10 streams
 * as the GPU engine (keyed by iteration, determinant index, attempt, purpose),
 * not from HANDE's dSFMT; stream-level parity with HANDE itself is therefore
 * unpinned, and whole runs are compared with the reference statistically.
 */
#ifndef HANDE_ORACLE_H
#define HANDE_ORACLE_H

#include <stdint.h>
#include "../include/hande_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_ctx oracle_ctx;

oracle_ctx *oracle_create(const hgpu_config *cfg, const hgpu_system *sys);
void oracle_destroy(oracle_ctx *c);
int oracle_initial_distribution(oracle_ctx *c);
int oracle_set_walkers(oracle_ctx *c, const int64_t *states, const int64_t *pops, const double *dat,
                       int64_t n);
int64_t oracle_get_walkers(oracle_ctx *c, int64_t *states, int64_t *pops, double *dat, int64_t cap);
int oracle_run_cycles(oracle_ctx *c, int32_t ncycles);
int oracle_end_report(oracle_ctx *c, hgpu_report *out);
int oracle_get_state(oracle_ctx *c, hgpu_state *out);
int oracle_set_state(oracle_ctx *c, const hgpu_state *in);
int oracle_eval_excitations(oracle_ctx *c, const int64_t *parents, const int64_t *parent_pops, int64_t n,
                            int64_t iteration, int32_t *orbs, double *pgen, double *hmatel,
                            int32_t *allowed, int64_t *nspawn);
int oracle_annihilate_fixed(oracle_ctx *c, const int64_t *sdata, int64_t n, int64_t iteration);
/* <D1|H|D2> (get_hmatel_hub_k / get_hmatel_mol) and <D|H|D> (sc0_ptr). */
double oracle_hmatel(oracle_ctx *c, const int64_t *f1, const int64_t *f2);
double oracle_sc0(oracle_ctx *c, const int64_t *f);
/* pgen of an explicit excitation (calc_pgen_* of the configured generator) */
double oracle_pgen(oracle_ctx *c, const int64_t *f, const int32_t *orbs);
/* pattempt_parallel of the spin-resolved generators (negative for the others). */
double oracle_pattempt_parallel(oracle_ctx *c);
/* pattempt_single and pattempt_double after init_excit_gen (src/qmc.F90:951-972). */
void oracle_pattempt(oracle_ctx *c, double *out);
/* The deterministic space of a semi-stochastic calculation (main-list order):
 * copied into dets when n is large enough; returns its size (0 before it is built). */
int64_t oracle_determ_space(oracle_ctx *c, int64_t *dets, int64_t n);
/* Replica 2-RDM (density_matrices): copies the current report's RDM
 * ([pair][pair], pairs p < q in tri_ind_distinct order) into out when n is
 * large enough and returns its element count (0 when not enabled); its
 * calc_rdm_energy; and, for tests, the diagonal contribution of the current
 * main list (update_rdm_from_spawns without spawns). */
int64_t oracle_rdm(oracle_ctx *c, double *out, int64_t n);
void oracle_rdm_energy(oracle_ctx *c, double *energy, double *trace);
void oracle_rdm_from_list(oracle_ctx *c);
/* Counters of the last cycles (spawn attempts etc.). */
int64_t oracle_total_attempts(oracle_ctx *c);
/* One calculation hash-partitioned over nthreads ranks (threads), as HANDE
 * runs it over MPI ranks: determinants owned by modulo(MurmurHash2, ranks),
 * spawned entries exchanged once per cycle, estimators summed per report.
 * Used to time the reference algorithm on all host cores. */
typedef struct oracle_par oracle_par;
oracle_par *oracle_par_create(const hgpu_config *cfg, const hgpu_system *sys, int nthreads);
void oracle_par_destroy(oracle_par *p);
int oracle_par_initial_distribution(oracle_par *p);
int oracle_par_begin_report(oracle_par *p);
int oracle_par_run_cycles(oracle_par *p, int32_t ncycles);
int oracle_par_end_report(oracle_par *p, hgpu_report *out);
int oracle_par_snapshot(oracle_par *p, int restore);
int oracle_par_set_state(oracle_par *p, const hgpu_state *in);
int oracle_par_get_state(oracle_par *p, hgpu_state *out);
int64_t oracle_par_total_attempts(oracle_par *p);
int64_t oracle_par_get_walkers(oracle_par *p, int64_t *states, int64_t *pops, double *dat, int64_t cap);
/* Philox4x32-10 uniform, for cross-checking the device generator. */
double oracle_uniform(uint64_t seed, uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, int which);

#ifdef __cplusplus
}
#endif

#endif
