/*
 * hande_gpu.h -- C ABI of the GB300 FCIQMC walker-propagation engine.
 *
 * The engine replaces the body of one FCIQMC Monte Carlo cycle of HANDE
 * (src/fciqmc.f90:307-399: init_mc_cycle, the loop over occupied
 * determinants with spawning and death, direct_annihilation, end_mc_cycle) and
 * the estimator/shift part of end_report_loop (src/qmc_common.F90:1082-1166 ->
 * src/energy_evaluation.F90:126-711) with kernels that run on one GPU, on
 * walker lists that stay resident in device memory between calls.
 *
 * Every entry point is extern "C", takes plain C scalars, pointers and POD
 * structs and returns an int status (HGPU_OK == 0), so the header can be bound
 * from Fortran with ISO_C_BINDING (bind(c) interfaces) as well as from C, C++
 * and Python ctypes.  No entry point aborts, traps or throws across the ABI.
 *
 * Conventions shared with HANDE's data model (src/qmc_data.f90:615-682,
 * lib/local/const.F90:25-56 with DET_SIZE=64, POP_SIZE=64):
 *   - a determinant is nwords = ceil(nbasis/64) int64 words; spin orbital p
 *     (0-based; HANDE orbital p+1) is bit p%64 of word p/64; even p are alpha
 *     (Ms=+1), odd p beta (src/basis_types.f90:134-170);
 *   - determinants are ordered by unsigned comparison with the LAST word most
 *     significant, ascending (src/bit_utils.F90:452-478, src/search.f90:47);
 *   - populations are int64 fixed point with pop_real_factor = 2^31 for real
 *     amplitudes and 1 otherwise (src/particle_t_utils.f90:53-82);
 *   - dat(1) of a walker is K_ii = <D_i|H|D_i> - E_HF (src/annihilation.f90:855).
 * Arrays passed across the ABI use HANDE's column-major layout: states(nwords, n)
 * i.e. the words of one determinant are contiguous, pops(nspaces, n).
 */
#ifndef HANDE_GPU_H
#define HANDE_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HGPU_MAX_WORDS 2   /* up to 128 spin orbitals */
#define HGPU_MAX_SPACES 2  /* nspaces: 1, or 2 with replica_tricks */

/* Status codes. */
enum {
    HGPU_OK = 0,
    HGPU_ERR_INVALID = 1,         /* invalid argument or configuration */
    HGPU_ERR_OOM = 2,             /* device allocation failed */
    HGPU_ERR_SPAWN_OVERFLOW = 3,  /* spawned list full (spawn%error, src/spawning.F90:938) */
    HGPU_ERR_MAIN_OVERFLOW = 4,   /* main list full (psip_list%error, src/annihilation.f90:750) */
    HGPU_ERR_TIMEOUT = 5,         /* a bounded device wait gave up */
    HGPU_ERR_CUDA = 6,            /* CUDA runtime error */
    HGPU_ERR_NO_DEVICE = 7,       /* no usable CUDA device */
    HGPU_ERR_UNSUPPORTED = 8      /* option outside what this build implements */
};

/* Error flags reported per report (bit mask). */
#define HGPU_FLAG_SPAWN_OVERFLOW 1
#define HGPU_FLAG_MAIN_OVERFLOW 2
#define HGPU_FLAG_TIMEOUT 4   /* a bounded device wait gave up (results of that cycle invalid) */
#define HGPU_FLAG_INTERNAL 8  /* an internal consistency check failed (results of that cycle invalid) */
#define HGPU_FLAG_BAD_DET 16  /* a spawned determinant has the wrong number of alpha or beta electrons
                                 (results of that cycle invalid) */

/* System kinds (sys%system in src/system.f90). */
enum { HGPU_SYS_HUB_K = 1, HGPU_SYS_READ_IN = 2 };

/* Excitation generators: same numbering as the excit_gen enum of
 * src/qmc_data.f90:31-68 (4 power_pitzer is not provided: HANDE itself refuses
 * it for read_in systems, src/check_input.F90:222-226). */
enum {
    HGPU_EXCIT_GEN_RENORM = 0,
    HGPU_EXCIT_GEN_RENORM_SPIN = 1,
    HGPU_EXCIT_GEN_NO_RENORM = 2,
    HGPU_EXCIT_GEN_NO_RENORM_SPIN = 3,
    HGPU_EXCIT_GEN_POWER_PITZER_OCC = 5,       /* 'uniform_power_pitzer' */
    HGPU_EXCIT_GEN_POWER_PITZER_OCC_IJ = 6,    /* 'heat_bath_power_pitzer' */
    HGPU_EXCIT_GEN_POWER_PITZER_ORDERN = 7,    /* 'heat_bath_power_pitzer_ref' */
    HGPU_EXCIT_GEN_CAUCHY_SCHWARZ_OCC = 8,     /* 'uniform_cauchy_schwarz' */
    HGPU_EXCIT_GEN_CAUCHY_SCHWARZ_OCC_IJ = 9,  /* 'heat_bath_cauchy_schwarz' */
    HGPU_EXCIT_GEN_HEAT_BATH = 10,
    HGPU_EXCIT_GEN_HEAT_BATH_UNIFORM = 11,
    HGPU_EXCIT_GEN_HEAT_BATH_SINGLE = 12
};

/* Arithmetic of the spawning step. */
enum {
    HGPU_PREC_FP64 = 0,   /* everything in FP64 (the reference's real(p) = real64) */
    HGPU_PREC_MIXED = 1   /* FP32 off-diagonal H_ij and p_gen; FP64 K_ii, shift, estimators */
};

/* The system, as HANDE holds it after init_system / read_in_integrals.  All
 * pointers are read during hgpu_create only (copied to device memory). */
typedef struct hgpu_system {
    int32_t kind;              /* HGPU_SYS_* */
    int32_t nbasis;            /* number of spin orbitals (sys%basis%nbasis) */
    int32_t nel, nalpha, nbeta;
    int32_t nwords;            /* ceil(nbasis/64) (sys%basis%tot_string_len) */
    const int32_t *orb_sym;    /* [nbasis] basis_fns(p+1)%sym: k-point index (hub_k) or irrep */
    const int32_t *orb_ms;     /* [nbasis] basis_fns(p+1)%ms: +1 or -1 */
    const double *sp_eigv;     /* [nbasis] single-particle eigenvalues */
    /* Hubbard model in momentum space (src/momentum_symmetry.f90:17-80). */
    int32_t nkpoints;          /* sys%nsym = nbasis/2 */
    const int32_t *sym_table;  /* [nkpoints*nkpoints] k_i+k_j, 0-based, row-major */
    const int32_t *inv_sym;    /* [nkpoints] -k_i, 0-based */
    double coulomb_k;          /* U/nsites (src/system.f90:578) */
    /* Molecular systems read from an FCIDUMP (src/read_in.F90, RHF, no Lz). */
    int32_t norb;              /* spatial orbitals M */
    int32_t nsym_pg;           /* number of irreps (power of two); cross product = XOR */
    const double *h1;          /* [norb*norb] one-body integrals, row-major, symmetric */
    const double *v2;          /* packed (ia|jb), index tri(tri(i,a),tri(j,b)); npair=M(M+1)/2 */
    int64_t nv2;               /* npair*(npair+1)/2 */
    double ecore;
    const int32_t *nbasis_sym_spin;    /* [2*nsym_pg] index ims*nsym_pg+sym; ims 0=beta 1=alpha */
    int32_t max_sym_spin;              /* max of nbasis_sym_spin */
    const int32_t *sym_spin_basis_fns; /* [nsym_pg*2*max_sym_spin] index (sym*2+ims)*max+k */
} hgpu_system;

/* Calculation options: the scalar fields of qmc_in_t / fciqmc_in_t
 * (src/qmc_data.f90:121-260) that the FCIQMC cycle uses. */
typedef struct hgpu_config {
    double tau;
    double shift_damping;          /* qs%shift_damping, default 0.05 */
    double initial_shift;
    double vary_shift_from;
    double target_particles;
    double initiator_pop;          /* initiator_threshold, default 3 */
    double spawn_cutoff;           /* in walker units (0.01 default) */
    double pattempt_single;        /* < 0: HANDE's default for the system */
    double pattempt_double;
    double D0_population;          /* init_pop */
    int32_t vary_shift_from_proje;
    int32_t excit_gen;             /* HGPU_EXCIT_GEN_* */
    int32_t real_amplitudes;
    int32_t initiator_approx;
    int32_t nspaces;               /* 1, or 2 for replica_tricks */
    int32_t ncycles;               /* mc_cycles per report */
    int32_t precision;             /* HGPU_PREC_* */
    int32_t quadrature_initiator;  /* fciqmc_in%quadrature_initiator (HANDE's default: 1): with two
                                      spaces the pair (N_1, N_2) of a determinant is an initiator in
                                      both iff N_1^2 + N_2^2 > initiator_pop^2 (set_parent_flag,
                                      src/ifciqmc.f90:14-57); 0: each space on its own */
    int64_t seed;                  /* rng_seed */
    int64_t walker_length;         /* main-list capacity; < 0 means MB (state_size) */
    int64_t spawned_walker_length; /* spawned-list capacity; < 0 means MB */
    uint64_t ref_det[HGPU_MAX_WORDS]; /* reference determinant f0 */
    double pattempt_parallel;      /* renorm_spin / no_renorm_spin: probability that a double
                                      excitation moves two electrons of parallel spin
                                      (choose_ij_spin_mol, src/excit_gen_mol.f90:684-783); < 0: the
                                      |H| ratio of find_parallel_spin_prob_mol
                                      (src/qmc_common.F90:265-378); > 0 with other generators is
                                      refused, as check_input does (src/check_input.F90:212-218) */
    int32_t density_matrices;      /* fciqmc_in%density_matrices: replica sampling of the 2-RDM
                                      (src/replica_rdm.F90); needs nspaces = 2, molecular systems */
    int32_t density_matrix_report; /* fciqmc_in%density_matrix_report: accumulate from the first
                                      report after this one in which every shift varies */
    double power_pitzer_min_weight;  /* qmc_in%power_pitzer_min_weight (HANDE's default 0.01):
                                        floor, as a share of the mean, of the weights of
                                        heat_bath_power_pitzer_ref's i, j and single tables
                                        (check_min_weight_ratio); must lie in [0, 1] */
    /* semi_stoch_in_t (src/qmc_data.f90:305-338) */
    int32_t semi_stoch_space;       /* space_type: 0 none, 1 'high' (the most populated
                                       determinants when the space is built), 4 'ci' (every
                                       determinant of the reference's spin and symmetry within
                                       semi_stoch_ci_level excitations of it; molecular systems) */
    int32_t semi_stoch_size;        /* target_size of a 'high' space */
    int64_t semi_stoch_start_iter;  /* start_iteration: the space is built at the start of
                                       this iteration (HANDE's default 1) */
    int64_t semi_stoch_shift_iter;  /* shift_start_iteration: built this many iterations after
                                       every shift varies (-1: not used) */
    int32_t semi_stoch_ci_level;    /* ci_space%ex_level of a 'ci' space */
    int32_t semi_stoch_combined;    /* 0: separate annihilation (HANDE's default: the projected
                                       amplitudes added to the main list); 1: combined
                                       (separate_annihilation = false: they join the spawned list
                                       as spawns from initiators, determ_proj_combined_annihil,
                                       src/semi_stoch.F90:897-975) */
    double shift_harmonic_forcing;  /* qs%shift_harmonic_forcing, the restoring factor zeta of the
                                       harmonic population control (update_shift,
                                       src/energy_evaluation.F90:659-711): every shift update also
                                       subtracts zeta ln(N_w / target_particles) / (tau A) when
                                       target_particles > 0; 0 gives the original dynamics */
    int32_t target_reference;       /* qmc_in%target_reference (the reference_target option): a
                                       shift starts to vary when its space's reference population
                                       N_0, not its total population, exceeds target_particles
                                       (communicated_energy_estimators,
                                       src/energy_evaluation.F90:638-650) */
    int32_t reserved0;
} hgpu_config;

/* One report line: the columns of write_qmc_report (src/qmc_io.f90:23-136). */
typedef struct hgpu_report {
    int64_t iteration;                       /* cycles completed so far */
    double shift[HGPU_MAX_SPACES];
    double proj_energy[HGPU_MAX_SPACES];     /* \sum H_0j N_j, averaged over the report */
    double D0_population[HGPU_MAX_SPACES];   /* N_0, averaged over the report */
    double nparticles[HGPU_MAX_SPACES];      /* # H psips at the end of the report */
    int32_t vary_shift[HGPU_MAX_SPACES];
    int64_t nstates;                         /* # states */
    int64_t nspawn_events;                   /* # spawn_events (last cycle) */
    double rspawn;                           /* R_spawn, averaged over cycles */
    int64_t nattempts;                       /* spawn attempts in the report (decide_nattempts sums) */
    int64_t nspawned;                        /* spawned entries in the report */
    int32_t error_flags;                     /* HGPU_FLAG_* */
    int32_t reserved0;
    double device_ms;                        /* device time of the report's cycles */
    double rdm_energy;                       /* RDM energy numerator of the report (calc_rdm_energy) */
    double rdm_trace;                        /* trace of the report's 2-RDM */
    /* bloom_stats_t (src/bloom_handler.F90:26-71, accumulate_bloom_stats :104):
     * spawning events that created at least 3 particles (the fixed-n threshold of
     * FCIQMC, src/fciqmc.f90:214) */
    int64_t nblooms;                         /* nblooms_curr: blooms in the report */
    double tot_bloom;                        /* tot_bloom_curr: particles created by them */
    double max_bloom;                        /* max_bloom: largest bloom of the calculation so far */
} hgpu_report;

typedef struct hgpu_handle hgpu_handle;

/* Library version (major*10000 + minor*100 + patch). */
int32_t hgpu_version(void);

/* Human-readable text for a status code. */
const char *hgpu_error_string(int32_t status);

/* Number of CUDA devices visible; 0 when no driver/device is present. */
int32_t hgpu_device_count(void);

/* Create an engine on the current CUDA device: copies the system to device
 * memory and allocates the main list, spawned list and scratch sized from
 * walker_length / spawned_walker_length.  Replaces init_qmc's allocation part
 * (src/qmc.F90:10-215, init_spawn_store :1418). */
int32_t hgpu_create(const hgpu_config *cfg, const hgpu_system *sys, hgpu_handle **out);

int32_t hgpu_destroy(hgpu_handle *h);

/* Put D0_population walkers on the reference determinant: initial_distribution
 * (src/qmc.F90:1507-1560); also sets the shift to initial_shift. */
int32_t hgpu_initial_distribution(hgpu_handle *h);

/* Replace the walker list.  states is (nwords, n) column-major, pops is
 * (nspaces, n) in encoded fixed point; dat may be NULL (K_ii is then
 * evaluated by slater_condon0).  The list must be sorted and unique. */
int32_t hgpu_upload_walkers(hgpu_handle *h, const int64_t *states, const int64_t *pops,
                            const double *dat, int64_t n);

/* Copy the walker list to the host.  *n_out receives the number of states;
 * nothing is written when capacity < *n_out (status HGPU_ERR_INVALID). */
int32_t hgpu_download_walkers(hgpu_handle *h, int64_t *states, int64_t *pops, double *dat,
                              int64_t capacity, int64_t *n_out);

/* The replica 2-RDM of the current report (density_matrices; the RDM array of
 * src/fciqmc.f90:134, rdm(p,q,r,s) in physical notation): rdm[row * npairs +
 * col] with npairs = nbasis (nbasis - 1) / 2, rows and columns the pairs
 * p < q of 0-based spin orbitals in tri_ind_distinct order (index q (q-1)/2 + p),
 * not normalised.  *n_out receives npairs^2 (0 without an RDM); rdm = NULL only
 * queries that size, and nothing is written when capacity is smaller
 * (HGPU_ERR_INVALID). */
int32_t hgpu_rdm_download(hgpu_handle *h, double *rdm, int64_t capacity, int64_t *n_out);

/* Run ncycles Monte Carlo cycles (src/fciqmc.f90:293-413) on the device;
 * estimators accumulate until hgpu_end_report. */
int32_t hgpu_run_cycles(hgpu_handle *h, int32_t ncycles);

/* Close a report loop: average the estimators over the cycles run since the
 * last call, update the shift and vary_shift (communicated_energy_estimators,
 * src/energy_evaluation.F90:425-657; update_shift :659-711). */
int32_t hgpu_end_report(hgpu_handle *h, hgpu_report *out);

/* Run one whole report (ncycles from the config, then hgpu_end_report). */
int32_t hgpu_run_report(hgpu_handle *h, hgpu_report *out);

/* Scalars of the qmc_state that a checkpoint needs. */
typedef struct hgpu_state {
    int64_t iteration;
    double shift[HGPU_MAX_SPACES];
    int32_t vary_shift[HGPU_MAX_SPACES];
    double nparticles_old[HGPU_MAX_SPACES];  /* N_w at the end of the last report */
    double tau;
    int64_t seed;
} hgpu_state;

int32_t hgpu_get_state(hgpu_handle *h, hgpu_state *out);
int32_t hgpu_set_state(hgpu_handle *h, const hgpu_state *in);

/* Write / read a binary checkpoint of the walker list and hgpu_state (the
 * logical fields of HANDE's restart file, src/restart_hdf5.F90:40-100, with
 * the counter-based RNG's (seed, iteration) in place of the dSFMT state). */
int32_t hgpu_checkpoint(hgpu_handle *h, const char *path);
int32_t hgpu_restore(hgpu_handle *h, const char *path);

/* ---- Parity entry points (fixed inputs, results returned to the host) ---- */

/* For n parent determinants (nwords each), draw one excitation with the
 * generator of the configuration, using RNG stream (iteration, parent index
 * i, attempt, space 0): gen_excit_ptr%full / %init+%finalise
 * (src/proc_pointers.f90:279-309).  Outputs per parent: from/to spin
 * orbitals (4 x int32, -1 when unused), p_gen, H_ij (signed), allowed flag,
 * and the encoded spawned population of the attempt (attempt_to_spawn,
 * src/spawning.F90:711) given parent_pops[i]. */
int32_t hgpu_eval_excitations(hgpu_handle *h, const int64_t *parents, const int64_t *parent_pops,
                              int64_t n, int64_t iteration, int32_t *orbs, double *pgen,
                              double *hmatel, int32_t *allowed, int64_t *nspawn);

/* Annihilate a fixed spawned list into the resident main list exactly as
 * direct_annihilation does (src/annihilation.f90:9-214): sort, self-annihilate
 * (src/spawn_data.F90:859/:937), annihilate_main_list[_initiator] (:294/:372),
 * remove_unoccupied_dets (:537), round_low_population_spawns (:600) and
 * insert_new_walkers (:677).  sdata is (nwords + nspaces + 1, n) column-major
 * (det words, pops, flag).  iteration keys the stochastic rounding. */
int32_t hgpu_annihilate_fixed(hgpu_handle *h, const int64_t *sdata, int64_t n, int64_t iteration);

/* K_ii = slater_condon0(D_i) - H00 for n determinants (sc0_ptr). */
int32_t hgpu_eval_diagonal(hgpu_handle *h, const int64_t *dets, int64_t n, double *kii);

/* Save (restore = 0) or restore (restore = 1) the walker list and the
 * population counters in device memory.  A benchmark or a caller that
 * replays cycles from one walker distribution restores it before each cycle
 * without a host round trip; the iteration counter keeps advancing, so every
 * replay draws fresh random numbers.  (No counterpart in the reference; its
 * nearest relative is reading a restart file, src/restart_hdf5.F90:539.) */
int32_t hgpu_snapshot(hgpu_handle *h, int32_t restore);

/* Self-annihilation of a spawned list with no device allocation by the
 * library.  For callers that cannot let a library allocate device memory: a
 * host program whose pool allocator owns all device memory, or a caller that
 * must not allocate on its critical path (cudaMalloc/cudaFree can synchronise
 * the device).  No counterpart in the reference.  The operation: sort the
 * entries by determinant (unsigned, last word most significant), add the
 * populations of equal determinants, drop the determinants whose populations
 * all cancel.
 *
 * d_sdata: device array (nwords + nspaces + 1, n) column-major, as for
 * hgpu_annihilate_fixed (the flag word is ignored); d_out: device array with
 * room for (nwords + nspaces, n) int64 -- receives the distinct determinants
 * in ascending order with their summed populations, entries whose populations
 * all cancel removed; *n_out (host): number of entries written.  stream: a
 * cudaStream_t, or NULL for the default stream; the call returns when the
 * work is done.
 *
 * Limits: n <= HGPU_NOALLOC_MAX_ENTRIES; larger lists are rejected with
 * HGPU_ERR_INVALID and *n_out = -HGPU_NOALLOC_MAX_ENTRIES.  The working space
 * is one fixed array (about 5 MB) inside the library, held on every GPU that
 * loads the library until the process exits.  The first call on a device looks
 * up that array's device address, so make it with that device current; the
 * address is kept for the life of the process, so a cudaDeviceReset between
 * calls (which destroys the context the address belongs to) is not supported.
 * Every call uses the same array: calls that overlap on the GPU (e.g. on two
 * streams or from two host threads) race; order them. */
#define HGPU_NOALLOC_MAX_ENTRIES 65536
int32_t hgpu_self_annihilate_noalloc(const int64_t *d_sdata, int64_t n, int32_t nwords, int32_t nspaces,
                                     int64_t *d_out, int64_t *n_out, void *stream);

/* Run one cycle with device timestamps between its phases (the role of
 * HANDE's per-section timing report, parallel_timing_t in
 * lib/local/parallel.F90:80-88).  phase_ms[0..6]: prep (E_proj, nattempts,
 * death), attempt scan, spawning, sort, self-annihilation, merge, end of
 * cycle.  counts[0..7] (may be NULL): N before, attempts, spawned, unique
 * spawned, N after, kernel launches per cycle, radix passes, bytes the radix
 * passes read and write per spawned entry (all passes together). */
int32_t hgpu_profile_cycle(hgpu_handle *h, double *phase_ms, int32_t nphase, int64_t *counts);

/* Launch shape of a handle's kernels (no counterpart in the reference, which
 * runs on CPU cores).  The results do not depend on it -- every count, sum and
 * random stream of a cycle is independent of how the work is split -- only the
 * speed does, so a caller (or an autotuner over a batch of handles) may change
 * it between cycles.  hgpu_create picks it from the list capacities.
 *   spawn_chunk    attempts a warp of the spawning kernel claims at a time:
 *                  32 to 256, a multiple of 32 (small chunks balance small
 *                  calculations, large ones cut the claims of large ones)
 *   spawn_blocks   blocks of the spawning kernel, >= 1
 *   stream_blocks  blocks of the streaming kernels (parent pass, scans,
 *                  annihilation, RDM), 1 to 1024
 *   sort_blocks    blocks of the radix-sort passes, >= 1
 * hgpu_set_launch rejects values outside these ranges (HGPU_ERR_INVALID). */
typedef struct hgpu_launch {
    int32_t spawn_chunk;
    int32_t spawn_blocks;
    int32_t stream_blocks;
    int32_t sort_blocks;
} hgpu_launch;

int32_t hgpu_get_launch(hgpu_handle *h, hgpu_launch *out);
int32_t hgpu_set_launch(hgpu_handle *h, const hgpu_launch *in);

/* Batches: many independent calculations advanced together.  HANDE runs one
 * calculation per process; a batch groups already-created handles (different
 * systems, sizes, seeds, replicas) on one device and advances all of them by
 * a cycle with a single CUDA graph launch, each handle's cycle a branch of the
 * graph, so small calculations fill the GPU together.  The handles stay owned
 * by the caller and must outlive the batch; hgpu_end_report and every other
 * per-handle call remain valid between batch calls.
 *
 * hgpu_batch_create: n >= 1 distinct handles on the current device.
 * hgpu_batch_run_cycles: ncycles cycles of every handle (as hgpu_run_cycles
 *   on each); handles must all be at the same buffer parity, which they are
 *   when they have run the same number of cycles since their list was set.
 *   Returns the first non-OK status of any handle (overflow flags), else OK.
 * hgpu_batch_destroy: frees the batch's graphs, not the handles. */
typedef struct hgpu_batch hgpu_batch;
int32_t hgpu_batch_create(hgpu_handle *const *handles, int32_t n, hgpu_batch **out);
int32_t hgpu_batch_run_cycles(hgpu_batch *b, int32_t ncycles);
int32_t hgpu_batch_destroy(hgpu_batch *b);

#ifdef __cplusplus
}
#endif

#endif /* HANDE_GPU_H */
