// hgpu_kernels.cuh -- device state and kernel launchers of one FCIQMC cycle.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "hgpu_device.cuh"

namespace hgpu {

constexpr int kBlock = 256;      // threads per block of the streaming kernels
// Largest chunk of attempts a warp claims from the spawning kernel's work
// counter (its queue size); the chunk of a handle (DevBuffers::spawn_chunk) is
// a multiple of 32 up to it.
constexpr int kSpawnChunk = 8 * 32;
// Generator kind of the spawning kernels (a template parameter, so that each
// kernel holds the code of one generator): HGPU_SYS_HUB_K, HGPU_SYS_READ_IN
// (molecular, uniform renorm generator) or one of the kinds below.
constexpr int kKindHeatBath = 3;         // molecular, heat_bath
constexpr int kKindReadInNoRenorm = 4;   // molecular, uniform no_renorm generator
constexpr int kKindHeatBathUniform = 5;  // molecular, heat_bath_uniform
constexpr int kKindPowerPitzerOcc = 6;   // molecular, uniform_ / heat_bath_ power_pitzer, cauchy_schwarz (FP64)
constexpr int kKindPowerPitzerRef = 7;   // molecular, heat_bath_power_pitzer_ref (FP64)
// pinfo bit of a main-list entry in the deterministic space (bits 0-1: sign of
// each space, 2-3: not an initiator in each space)
constexpr uint8_t kDetermBit = 0x80;
// Radix sort of the spawned list (hgpu_sort.cuh): 8-bit digits, at most
// kMaxPasses passes, tiles of kOSThreads x items keys of KW words each.
constexpr int kOSThreads = 256;  // one thread per digit value in the look-back
constexpr int kMaxPasses = 16;
template <typename K, int KW>
struct OSConf {
    // keys per thread (4 blocks of 256 fit an SM)
    static constexpr int items = sizeof(K) * KW <= 8 ? 12 : 6;
    static constexpr int tile = kOSThreads * items;
    static constexpr size_t smem = (size_t)tile * (sizeof(K) * KW + 4);  // staged keys + indices
};
constexpr int kRadixBits = 8;
constexpr int kRadix = 1 << kRadixBits;
constexpr int kSortItems = 8;    // keys per thread per radix tile
constexpr int kMaxBlocks = 1024; // upper bound of the fixed grid (partials arrays)
// Merged elements per annihilation tile (hgpu_annihilate.cu): 2048 for one-word
// determinants, 1024 for two-word ones, whose tiles take twice the shared
// memory per element; kAnnTileMin sizes the per-tile arrays.
template <int W>
constexpr int ann_tile() {
    return W == 1 ? 2048 : 1024;
}
constexpr int kAnnTileMin = 1024;
// Bloom threshold of FCIQMC in particles: init_bloom_stats_t's default with
// bloom_mode_fixedn (src/fciqmc.f90:214, src/bloom_handler.F90:37).
constexpr int64_t kBloomThreshold = 3;

// Per-cycle counters and per-report accumulators, resident in device memory so
// that a whole cycle runs without host synchronisation (and can be replayed
// as a CUDA graph).  Sizes of the variable-length lists live here.
struct DevState {
    int64_t n_main;        // N: occupied determinants
    int64_t n_spawn;       // S: spawned entries this cycle
    int64_t n_uniq;        // U: spawned determinants with a non-zero summed population
    int64_t n_attempts;    // A: spawning attempts this cycle
    int64_t n_merged_keep; // uint2 (kept main, kept total) after the annihilation
    int64_t n_slots;       // N * nspaces
    int64_t iter;          // current iteration (cycle number, 1-based)
    double shift[HGPU_MAX_SPACES];
    int64_t abs_pop[HGPU_MAX_SPACES];  // exact sum |pop| of the main list (encoded units)
    int64_t nattempts_cycle;           // nint(2 N_w) at the start of the cycle (rspawn)
    int32_t error_flags;
    int32_t pad;
    // report accumulators
    double acc_proj[HGPU_MAX_SPACES], acc_proj_c[HGPU_MAX_SPACES];
    double acc_d0[HGPU_MAX_SPACES], acc_d0_c[HGPU_MAX_SPACES];
    double acc_rspawn;
    int64_t acc_attempts, acc_spawned, last_nspawn_events;
    int32_t rep_cycles;
    int32_t pad2;
    uint64_t spawn_next;  // next unclaimed attempt chunk of the spawning kernel
    int64_t n_sq;         // singles queued for the singles kernel (may pass sq_cap: see k_spawn)
    int64_t n_spawn_stoch; // spawned entries from spawning attempts (the rest, with combined
                           // semi-stochastic annihilation, are the deterministic projection's)
    uint32_t os_ticket[16];  // next tile of each radix pass (hgpu_sort.cuh)
    uint32_t ann_ticket[2];  // next tile of each annihilation pass (hgpu_annihilate.cu)
    // replica 2-RDM (hgpu_rdm.cu)
    int32_t rdm_on;          // spawn_rdm active (set by the host at a report's start)
    int32_t pad4;
    int64_t n_rdm;           // RDM spawns of the cycle
    double rdm_energy, rdm_trace;  // calc_rdm_energy of the report
    // bloom_stats_t (src/bloom_handler.F90:26-71): spawning events of at least
    // kBloomThreshold particles -- their number and summed |amount| (encoded)
    // in the report, the largest |amount| of the calculation
    int64_t bloom_n, bloom_tot;
    uint64_t bloom_max;
};

// Device buffers of one engine (all allocated once, at create).
struct DevBuffers {
    // main list, double-buffered: states (nw per entry), pops (R per entry), K_ii
    uint64_t *dets[2];
    int64_t *pops[2];
    double *kii[2];
    int64_t cap;
    // per-parent work arrays (size cap)
    uint32_t *natt;     // attempts per (parent, space)
    int64_t *aoff;      // inclusive offsets of natt
    uint8_t *pinfo;     // per parent: bit s = sign(pop_s) < 0, bit 2+s = non-initiator in space s
    // spawned list (size scap)
    uint64_t *sdets;
    int64_t *spops;
    uint64_t *sflag;    // initiator bits | generation order << 2
    int64_t scap;
    // singles of the generators that draw the single/double choice first:
    // (slot, attempt in slot, stream position) queued by the spawning kernel
    // for the singles kernel (null for the other generators)
    uint4 *sq;
    int64_t sq_cap;
    // sort (hgpu_sort.cuh)
    uint64_t *skeys;    // ranks of the spawned determinants (when use_rank; 32-bit words when key32)
    uint64_t *keys[2];  // key_words per entry (32-bit words when key32)
    uint32_t *idx[2];
    uint32_t *ghist;    // [kMaxPasses][kRadix] digit counts
    uint32_t *gofs;     // [kMaxPasses][kRadix] global digit offsets
    uint64_t *lookback; // [tiles][kRadix] look-back status words
    uint32_t *os_epoch;  // look-back epoch of the current sort (kept out of DevState,
                         // which the host rewrites, so that an epoch is never reused)
    const uint64_t *binom;  // rank table [binom_rows][binom_cols] (hgpu_sort.cuh, det_rank)
    int use_rank;       // keys are ranks (1: one table load per electron, 2: two loads and a
                        // product, 3: the same with 128-bit products, two key words); 0: the
                        // keys are the determinant words
    int key32;          // the ranks fit 32 bits: 32-bit keys
    int key_words;
    int binom_rows, binom_cols;  // shape of the rank table
    int sort_na, sort_nb;        // electrons of each spin of every determinant
    int sort_few_from;          // first pass whose digits take at most 32 values
    int sort_few_values[16];    // number of digit values of each such pass
    int sort_grid;      // blocks of the radix passes
    int sort_packed;    // ranks sorted as packed records (hgpu_sort.cuh, P64 / P128): 0 no, else the
                        // words of the first record (1 or 2)
    int sort_key_bits;  // bits of the rank keys
    int sort_ibits;     // bits of the entry index in a packed record
    // annihilation (hgpu_annihilate.cuh)
    int64_t *msplit;       // per tile boundary: main index, spawned index, spawned index at the group boundary
    uint64_t *seg_status;  // per annihilation tile: look-back status word
    uint32_t *seg_epoch;   // look-back epoch of the annihilation (kept out of DevState)
    int splits_grid;       // blocks of k_ann_splits
    // replica 2-RDM (hgpu_rdm.cu; null unless density_matrices)
    double *rdm;            // [npairs][npairs], pairs p < q in tri_ind_distinct order
    int64_t npairs;
    uint64_t *rdm_schild;   // per RDM spawn: the child's words (size scap)
    uint32_t *rdm_sparent;  // per RDM spawn: the parent's index in the cycle's (old) main list
    int64_t *rdm_spops;     // per RDM spawn: amount
    uint8_t *rdm_sspace;    // per RDM spawn: space of the parent
    double *rdm_rows;       // [2][npairs]: per-row energy and diagonal of calc_rdm_energy
    uint32_t *rdm_hash;     // open-addressing table of the new main list (index per slot)
    int64_t rdm_hash_mask;  // table size - 1 (a power of two, at least 1.5 x cap)
    uint32_t rdm_hash_tagmask;  // entry bits above the list index: a tag from the hash's high word
    // the RDM diagonal runs on a second stream beside the RDM spawns (host
    // handles: a fork and a join event around it)
    cudaStream_t rdm_aux;
    cudaEvent_t rdm_fork, rdm_join;
    // semi-stochastic projection (hgpu_semi_stoch.cu): the deterministic
    // determinants in main-list order, the Hamiltonian by column j (rows i
    // ascending: H(D_i, D_j), diagonal K_jj), the populations of the
    // deterministic states at the start of the cycle ([nd][R], walker units)
    // and their main-list positions; nd = 0 until the space is built
    const uint64_t *ddets;
    const int64_t *dcol_ptr;
    const int32_t *dcol_i;
    const double *dcol_h;
    double *dvec;
    int64_t *dind;
    int64_t nd;
    int ss_combined;        // combined annihilation: the projection goes to the spawned list
    // scan scratch and per-block partials
    int64_t *scan_part;     // kMaxBlocks * 2
    double *part_d;         // kMaxBlocks * 4 (proj, d0 per space)
    int64_t *part_i;        // kMaxBlocks * 4 (abs pop per space, ndeath)
    DevState *state;
    DevSys *sys;
    int grid;               // blocks of the streaming kernels (at most kMaxBlocks)
    int spawn_grid;         // blocks of the spawning kernel
    int spawn_chunk;        // attempts a warp of the spawning kernel claims at a time (32..256, x32)
    int sort_passes;
    size_t fx_smem_bytes;  // exact-diagonal tables staged by the annihilation tiles (0: read
                           // through the L1 cache from global memory, for tables too large to
                           // stage without costing resident blocks)
    int nk;                 // hub_k: number of k-points (shared-memory tables)
};

// Events recorded between the phases of a cycle in profiling mode:
// 0 start, 1 after prep, 2 after attempt scan, 3 after spawn, 4 after sort,
// 5 after the merge-path cuts, 6 after the annihilation, 7 end.
constexpr int kNumMarks = 8;
struct PhaseMarks {
    cudaEvent_t ev[kNumMarks];
};

// One cycle, split in launchable phases.  cur = buffer index of the main list
// at the start of the cycle; the merged list is written to 1-cur.
void launch_cycle(const DevBuffers &b, int W, int R, int kind, int precision, int cur, cudaStream_t st,
                  const PhaseMarks *pm = nullptr);
int launches_per_cycle(const DevBuffers &b);
// Kernel attributes that depend on the system (dynamic shared memory); 0 on success.
int set_kernel_attributes(const DevBuffers &b);
void launch_annihilation(const DevBuffers &b, int W, int R, int kind, int cur, cudaStream_t st);
// Sort and annihilation of one cycle (hgpu_annihilate.cu), and the kernel
// attributes they need; 0 on success.
void launch_sort_annihilate(const DevBuffers &b, int W, int R, int cur, cudaStream_t st, const PhaseMarks *pm);
int set_annihilate_attributes(const DevBuffers &b);
// hgpu_semi_stoch.cu: the deterministic Hamiltonian by column (count, then fill
// at the offsets dcol_ptr), and each cycle's deterministic projection added to
// the main list
void launch_determ_columns(const DevBuffers &b, int W, int kind, bool fill, int64_t *counts, int32_t *col_i,
                           double *col_h, cudaStream_t st);
void launch_determ_project(const DevBuffers &b, int R, int cur, cudaStream_t st);
void launch_eval_excitations(const DevBuffers &b, int W, int kind, int precision, const uint64_t *parents,
                             const int64_t *parent_pops, int64_t n, int64_t iteration, int32_t *orbs, double *pgen,
                             double *hmatel, int32_t *allowed, int64_t *nspawn, cudaStream_t st);
void launch_eval_diagonal(const DevBuffers &b, int W, const uint64_t *dets, int64_t n, double *kii, cudaStream_t st);
void launch_load_fixed_spawns(const DevBuffers &b, int W, int R, const int64_t *sdata, int64_t n, cudaStream_t st);
void launch_abs_pop(const DevBuffers &b, int R, int cur, cudaStream_t st);
// Replica 2-RDM (hgpu_rdm.cu): the cycle's RDM spawns and diagonal into b.rdm
// (main list in buffer cur), calc_rdm_energy into DevState, kernel attributes.
void launch_rdm_cycle(const DevBuffers &b, int W, int R, int cur, cudaStream_t st);
// The spawning kernel of molecular systems that also records the RDM spawns
// (hgpu_spawn_rdm.cu); sm = its dynamic shared memory.
void launch_spawn_rdm(const DevBuffers &b, int W, int R, int kind, int precision, int cur, size_t sm,
                      cudaStream_t st);
void launch_rdm_energy(const DevBuffers &b, int W, cudaStream_t st);
int set_rdm_attributes();

}  // namespace hgpu
