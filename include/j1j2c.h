/*
 * libj1j2cuda — GB300 (sm_103a) Monte Carlo engine for the hot path of sim/J1J2_6tv.f90
 * (ShadowQFT/J1J2-public): single-spin Metropolis sweeps of the L x L x H J1-J2-Jperp model with
 * the random field on the nematic variable, the parallel-tempering (PT) swap, the observable
 * reductions and the per-slot running sums.  All disorder configurations ("confs") and all
 * replicas of their temperature ladders stay resident on one GPU.
 *
 * C ABI: plain pointers and sizes, int status (0 = OK, negative = error, text in
 * j1j2c_last_error).  Host arrays are caller-owned and are copied during the call; no pointer is
 * kept after a call returns.  Site order of every per-site array is the reference's
 * site = ix + L*iy + L*L*iz (J:539).  Replica, slot and pair indices are 0-based (the Fortran
 * binding adds 1).  Calls are synchronous at return unless stated otherwise.
 *
 * Each entry point names the reference code it replaces ("J:" = sim/J1J2_6tv.f90,
 * "CR:" = sim/corr_rand_3d.f90).
 */
#ifndef J1J2C_H
#define J1J2C_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes (argument checks mirror Validate_run_options, J:841-925) */
#define J1J2C_OK 0
#define J1J2C_EINVAL -1   /* bad argument: odd L or H, NREPLICA != ladder size, bad enum ...    */
#define J1J2C_ECUDA -2    /* CUDA runtime error (text in j1j2c_last_error)                      */
#define J1J2C_ETIMEOUT -3 /* a bounded device wait expired                                      */
#define J1J2C_ENOMEM -4   /* device or host allocation failed                                   */
#define J1J2C_ESTATE -5   /* call order: e.g. run before every conf has disorder and a ladder  */

/* precision of the sweep (the swap, energies and running sums are FP64 in both forms) */
#define J1J2C_FP64_PLAIN 0   /* FP64 field and acceptance, bit-identical to the host replay      */
#define J1J2C_FP32_BATCHED 1 /* FP32 field and acceptance (ln u < -beta dE form)                 */

/* START / STRAXIS (J:62-63, Initialize_spin_array J:1179-1209) */
#define J1J2C_START_HOT 0 /* device Philox stream: s = +1 when u < 1/2                           */
#define J1J2C_START_FER 1
#define J1J2C_START_STR 2
#define J1J2C_AXIS_X 0 /* stripes run along x: s = (-1)^iy */
#define J1J2C_AXIS_Y 1 /* stripes run along y: s = (-1)^ix */

/* j1j2c_params.flags */
#define J1J2C_FLAG_NO_GRAPH 1u   /* launch kernels directly instead of replaying a CUDA graph     */
#define J1J2C_FLAG_PROFILE 2u    /* time every sweep launch with CUDA events (j1j2c_get_profile)  */
#define J1J2C_FLAG_GENERIC 4u    /* force the per-site kernel path (testing)                      */
#define J1J2C_FLAG_NO_FIXED 8u   /* skip the shape-specialised kernels (testing)                  */
#define J1J2C_FLAG_GLOBAL 16u    /* force the global-memory (one launch per colour) path (testing) */
#define J1J2C_FLAG_CLUSTER 64u   /* force the thread-block-cluster path, largest cluster that fits
                                    (testing; with J1J2C_FLAG_GENERIC one site per thread)        */
#define J1J2C_FLAG_WOLFF 32u     /* one Wolff cluster update at the start of every PT cycle       */
#define J1J2C_FLAG_WOLFF_SPLIT 1024u /* with J1J2C_FLAG_WOLFF and lattices in HBM (one launch per
                                        colour): the Wolff update and sweeps of the coldest quarter
                                        of the slots on one stream, those of the other slots on a
                                        second one; J1J2C_SPLIT="k1,k2,..." in the environment
                                        splits the slots at k1, k2, ... into up to eight ranges on
                                        as many streams (testing; else tuned)                     */
#define J1J2C_FLAG_STREAM 512u   /* the streaming form of the shape-specialised kernels: one CTA
                                    per SM through a range of lattices (testing; else tuned)      */
#define J1J2C_FLAG_WOLFF_BITS 2048u /* the Wolff growth reads bond activations decided beforehand
                                        for every lattice on every SM (testing; else tuned for the
                                        coldest slots of the split form)                          */
#define J1J2C_FLAG_PAIRS 4096u   /* the shape-specialised kernels with two replicas of one
                                    configuration per CTA, sharing the field copy (testing; else
                                    tuned)                                                        */
#define J1J2C_FLAG_MULTI 8192u   /* several lattice-shape groups (L = H = 16, 24, 32, 48): every
                                    group's sweeps in one persistent launch (testing; else tuned
                                    against one graph branch per group)                          */
#define J1J2C_FLAG_COOP 16384u   /* small batches: every colour phase, sweep and the observables of
                                    a cycle in one cooperative launch with grid barriers between
                                    the phases (testing; slower than one launch per phase,
                                    never chosen by the tuner)                                   */
#define J1J2C_FLAG_REPLICA 32768u /* small batches: the lattice replicated in every CTA of a
                                     thread-block cluster (the largest of 16, 8, 4, 2 CTAs that
                                     fits), every sweep and the observables of a cycle in one
                                     launch (testing; slower than one launch per phase, never
                                     chosen by the tuner)                                        */
#define J1J2C_FLAG_WOLFF_ASYNC 65536u /* one-CTA Wolff growths in the level-free form (a work
                                         queue instead of breadth-first levels; testing: no
                                         faster, never chosen by the tuner)                     */
#define J1J2C_FLAG_WOLFF_CS2 128u /* Wolff growth over 2 CTAs per lattice (testing; else tuned)    */
#define J1J2C_FLAG_WOLFF_CS4 256u /* Wolff growth over 4 CTAs per lattice (testing; else tuned);
                                     both flags: 2 CTAs for the coldest quarter of the slots, one
                                     for the rest                                                  */

/* Run parameters: the compile-time constants of J:43-96 that the hot path consumes. */
typedef struct {
    int32_t L, H;          /* lattice (both even: the 8-colour update needs it)                  */
    double J1h, J1v;       /* nearest-neighbour couplings along x and y (J1 +/- deltaJ1)        */
    double J2, J3;         /* diagonal and inter-layer couplings                                 */
    int32_t nconf;         /* disorder configurations resident in this context                  */
    int32_t nreplica;      /* PT ladder length per conf (NREPLICA = NTEMP); 1 = LOCAL sampler   */
    int32_t ptswapever;    /* sweeps per PT cycle (PTSWAPEVER)                                   */
    int32_t precision;     /* J1J2C_FP64_PLAIN or J1J2C_FP32_BATCHED                             */
    uint32_t seed;         /* Philox key word 0 (IRINIT)                                         */
    uint32_t conf_base;    /* Philox key word 1 of conf 0 (conf c uses conf_base + c)           */
    int32_t device;        /* CUDA device ordinal                                                */
    uint32_t flags;        /* J1J2C_FLAG_*                                                       */
    int32_t block_threads; /* 0 = autotuned; otherwise threads per CTA (multiple of 32, <=1024;
                              with lattices in HBM, one of the HBM kernel's sizes 128, 256,
                              512 where it has that shape)                                   */
} j1j2c_params;

/* Per (conf, slot) running sums of Pt_measurement_loop (J:1440-1513), in this order. */
typedef struct {
    double mag, absmag, mag2, mag4;
    double en, en2;
    double strx_abs, stry_abs, strx2, strx4, stry2, stry4;
    double str2, str4, absstr, nem;
    double nbar, nbarabs, nbar2, nbar4;
    double best_en, final_en;
    int64_t nmeasure;
} j1j2c_slot_sums;

/* Run description for the reference-format output files (the parameters Write_files prints,
 * J:43-96); strings are the reference's values, e.g. impmode "RAN", start "HOT", straxis "X",
 * samplermode "PT   ", updateorder "SEQ", tempprotocol "INDEP", ptstartmode "COMMON",
 * ptladdermode "LINEAR". */
typedef struct j1j2c_run_info {
    int32_t L, H;
    double J1, deltaJ1, J2, J3, phi, xi, pp;
    const char *impmode, *start, *straxis, *samplermode, *updateorder, *tempprotocol,
        *ptstartmode, *ptladdermode;
    int32_t nreplica, ptswapever, ptmeasindex, nconf, neq, nmess, irinit;
    double tladdermid, tladderfrac;
    int32_t bins;            /* BINS: > 0 writes the histogram file cfhs */
    int32_t write_strip;     /* WRITESTRIP: per-configuration stripe file cfxy */
    int32_t write_numflips;  /* WRITENUMFLIPS: per-site flip counts cfnu */
    int32_t write_phitable;  /* WRITEPHITABLE: random field table cfph */
} j1j2c_run_info;

/* Optional diagnostics of measured PT cycles (all off in a new context). */
typedef struct j1j2c_diagnostics {
    int32_t locnem_slot;  /* >= 0: per-site sums of s and of the local nematic term of the replica
                             at this slot (PTMEASINDEX - 1) after every measured cycle; -1: off */
    int32_t hist_bins;    /* > 0: per-slot energy histogram with this many bins (BINS); 0: off */
    int32_t trace_cycles; /* > 0: record {mag, en, strx, stry, nbar} of every slot and temp_of_rep
                             of every replica for the first trace_cycles measured cycles */
    int32_t flip_counts;  /* 1: per-site accepted flips per temperature slot; 0: off */
} j1j2c_diagnostics;

/* ---------------------------------------------------------------------------------------------
 * Context life cycle
 * ------------------------------------------------------------------------------------------- */

/* Allocates every device buffer for nconf x nreplica lattices.  Replaces the MPI set-up and the
 * per-rank arrays (J:115-207, Setup_mpi J:415-420, Setup_neighbor_table J:532-586). */
int j1j2c_create(void **ctx, const j1j2c_params *params);

/* Mixed lattice shapes in one context (one graph per PT cycle covers every group): group k
 * contributes groups[k].nconf confs of groups[k].L x L x H with groups[k].nreplica replicas;
 * confs are numbered across groups in order.  Couplings, ptswapever, precision, seed,
 * conf_base, device and flags are taken from groups[0]; block_threads is per group.  No
 * reference counterpart: the reference runs one lattice size per build (J:43-44). */
int j1j2c_create_multi(void **ctx, const j1j2c_params *groups, int32_t ngroups);

/* Lattice extents and ladder length of one conf (useful with j1j2c_create_multi). */
int j1j2c_conf_shape(void *ctx, int32_t conf, int32_t *L, int32_t *H, int32_t *nreplica);

/* Frees everything (J:401 MPI_FINALIZE's role for this context). */
void j1j2c_destroy(void *ctx);

/* Text of the last error on this context (or of the last failed create when ctx is NULL). */
const char *j1j2c_last_error(void *ctx);

/* Use a caller-provided cudaStream_t for all later work (NULL = the context's own stream). */
int j1j2c_set_stream(void *ctx, void *cuda_stream);

/* ---------------------------------------------------------------------------------------------
 * Inputs (replace the per-config set-up that feeds the hot path)
 * ------------------------------------------------------------------------------------------- */

/* Disorder of one conf: random field p (N doubles), occupancy (N int8, NULL = all occupied),
 * bond masks jh / jv (N int8, NULL = all bonds present).  Replaces the arrays filled by
 * Setup_vacancies (J:1111-1165) and Setup_phi_table (J:590-633) as the sweep reads them. */
int j1j2c_set_disorder(void *ctx, int32_t conf, const double *p, const int8_t *occu,
                       const int8_t *jh, const int8_t *jv);

/* Inverse temperatures of the ladder slots of one conf (NREPLICA doubles, slot 0 = TMIN);
 * conf < 0 sets every conf from nconf x NREPLICA doubles.  Replaces beta_ladder
 * (Setup_temperature_ladder J:928-962). */
int j1j2c_set_ladder(void *ctx, int32_t conf, const double *beta);

/* Initial spins of every replica of a conf, identity slot maps and zeroed swap counters.
 * spins == NULL generates START/STRAXIS (HOT from the device Philox stream); otherwise spins
 * holds NREPLICA x N int8 (+1/-1, replica-major).  Vacancies are stored as 0.  Must follow
 * j1j2c_set_disorder of the conf.  Replaces Initialize_pt_state (J:1218-1247) /
 * Initialize_spin_array (J:1179-1209). */
int j1j2c_init_spins(void *ctx, int32_t conf, int32_t start, int32_t axis, const int8_t *spins);

/* Zero the running sums, measurement counts and visit flags of one conf (conf < 0: all) and
 * reset best_en to +inf, as at the start of Pt_measurement_loop (J:1361-1389, J:1394-1395).
 * Swap counters run on across both loops, as cfg_ptswap_* do (reset by j1j2c_init_spins). */
int j1j2c_reset_measurements(void *ctx, int32_t conf);

/* Enable / disable the measurement diagnostics (replaces the WRITELOCNEM, WRITEHIST,
 * WRITEBINDTIME / trace and WRITENUMFLIPS bookkeeping of J:1009-1025, J:1397-1477,
 * J:1514-1523, J:1168-1177 and J:2575).  Every enabled diagnostic starts from zero.  Flip
 * counting runs the generic sweep kernels (the shape-specialised ones do not count) and is
 * charged 8 bytes of traffic per accepted flip; the others cost one small kernel or a few
 * stores per measured cycle.  The local nematic sums and the histogram restart with
 * j1j2c_reset_measurements (J:1388, J:1227-1230); flip counts restart with j1j2c_init_spins
 * (J:1231-1232); the trace is indexed by the measured-cycle count. */
int j1j2c_set_diagnostics(void *ctx, const j1j2c_diagnostics *diag);

/* ---------------------------------------------------------------------------------------------
 * Hot path
 * ------------------------------------------------------------------------------------------- */

/* ncycles PT cycles over every conf: PTSWAPEVER sweeps of every replica at its slot's beta, the
 * observable reduction of every replica, the alternating odd/even adjacent swap and (measure != 0)
 * the visit flags and per-slot running sums.  restart_swap_phase != 0 starts with pairs
 * (0,1),(2,3),... as both PT loops do (J:1266, J:1429).  Replaces Pt_equilibration_loop
 * (J:1250-1279) and the cycle loop of Pt_measurement_loop (J:1428-1532); with NREPLICA = 1 and
 * PTSWAPEVER = 1 it is the LOCAL Equilibration_loop / Measurement_loop (J:2122-2216). */
int j1j2c_run(void *ctx, int32_t ncycles, int32_t measure, int32_t restart_swap_phase);

/* The same cycles enqueued on the context's stream without waiting for them (j1j2c_run is this
 * followed by j1j2c_sync): the caller overlaps host work or queues further stream work behind
 * them.  Until j1j2c_sync returns, no other call may read or change the context's state. */
int j1j2c_enqueue(void *ctx, int32_t ncycles, int32_t measure, int32_t restart_swap_phase);

/* Waits for every enqueued cycle and reports as j1j2c_run does (J1J2C_ETIMEOUT when a bounded
 * device wait gave up, the context staying usable). */
int j1j2c_sync(void *ctx);

/* Drop-in for one call of Metro_sweep (J:2544-2608) on one lattice: nsweeps FP64 sweeps of
 * replica rep of conf at inverse temperature beta, Philox sweep counter starting at sweep_index.
 * On return mag/en/strx/stry (each may be NULL) hold the Measurement values (J:2807-2842) of the
 * new configuration; Fortran callers pass their curmag/curen/curstrx/curstry. */
int j1j2c_metro_sweep_fp64(void *ctx, int32_t conf, int32_t rep, double beta,
                           uint32_t sweep_index, int32_t nsweeps, double *mag, double *en,
                           double *strx, double *stry);

/* One Wolff cluster update of every lattice at its slot's beta: bonds with K s_i s_j > 0 are
 * activated with probability 1 - exp(-2 beta K s_i s_j) (K the per-bond coupling of
 * Compute_local_field, J:2498-2541) and the cluster of a Philox-chosen seed site is flipped.
 * By default one CTA per lattice grows the seed's cluster breadth-first; J1J2C_FLAG_NO_FIXED
 * selects shared-memory slab union-find labelling and J1J2C_FLAG_GENERIC per-site global
 * union-find labelling (scratch the context allocates on first use); all three flip the same
 * cluster.
 * The random stream is indexed by the PT cycle counter (a cycle with J1J2C_FLAG_WOLFF runs this
 * before its sweeps).  cluster_sizes (NULL or nconf x NREPLICA) receives the flipped sizes.
 * Replaces the Wolff update named in the reference's header (J:7), which it never implements. */
int j1j2c_wolff(void *ctx, int64_t *cluster_sizes);

/* Attempts per bond that the union-find labelling forms of the Wolff update (J1J2C_FLAG_NO_FIXED,
 * J1J2C_FLAG_GENERIC) make to merge two clusters before giving up (default 2^20, tries >= 0).
 * A labelling that gives up flips a cluster that may be incomplete, and the call that ran it
 * (j1j2c_wolff, or j1j2c_run with J1J2C_FLAG_WOLFF) returns J1J2C_ETIMEOUT; the error is then
 * cleared and the context stays usable.  For tests of that path (0 makes every activated bond
 * give up); no reference counterpart (the reference stops on errors, J:443-444). */
int j1j2c_set_retry_budget(void *ctx, int32_t tries);

/* Flipped-cluster sizes of the last Wolff update of one conf (NREPLICA; conf < 0: all). */
int j1j2c_get_cluster_sizes(void *ctx, int32_t conf, int64_t *out);

/* Deterministic replay audit of the FP32 form: nsweeps FP64 sweeps of every lattice at its slot's
 * beta, evaluating at every attempt the FP32 decision on the same configuration and uniform.
 * Adds to *attempts and *mismatches (FP32 decision != FP64 decision).  No reference
 * counterpart: it quantifies the FP32 form's deviation from the FP64 acceptance of J:2572-2604. */
int j1j2c_audit_fp32(void *ctx, int32_t nsweeps, int64_t *attempts, int64_t *mismatches);

/* ---------------------------------------------------------------------------------------------
 * Outputs
 * ------------------------------------------------------------------------------------------- */

/* Running sums of every slot of a conf (NREPLICA records; conf < 0: nconf x NREPLICA). */
int j1j2c_get_slot_sums(void *ctx, int32_t conf, j1j2c_slot_sums *out);

/* Swap attempts / accepts per adjacent pair (NREPLICA-1 each, may be NULL) and the number of
 * replicas that visited both ladder ends while measuring (cfg_ptswap_* and cfg_ptvisitboth,
 * J:1303-1338, J:1537). */
int j1j2c_get_pt_stats(void *ctx, int32_t conf, int64_t *attempts, int64_t *accepts,
                       int32_t *visited_both);

/* Slot maps rep_at_temp / temp_of_rep (NREPLICA each, 0-based; either may be NULL). */
int j1j2c_get_maps(void *ctx, int32_t conf, int32_t *rep_at_temp, int32_t *temp_of_rep);

/* Spins of one replica (N int8 in site order; vacancies read 0). */
int j1j2c_get_spins(void *ctx, int32_t conf, int32_t rep, int8_t *out);

/* Observables of every replica after the last cycle: NREPLICA x {mag, en, strx, stry, nbar}
 * (per occupied site; en includes the phi term, J:2835-2840; nbar as J:1028-1048);
 * conf < 0: every conf, nconf x NREPLICA x 5. */
int j1j2c_get_observables(void *ctx, int32_t conf, double *out);

/* Current diagnostics settings of the context. */
int j1j2c_get_diagnostics(void *ctx, j1j2c_diagnostics *out);

/* Occupied sites of one conf (N - nimp of its disorder; N before j1j2c_set_disorder). */
int j1j2c_get_occupied(void *ctx, int32_t conf, int32_t *nocc);

/* Per-site sums of the local nematic average of one conf (N doubles each, site order, either
 * may be NULL) and the number of cycles they hold: locspin_accum, locnem_accum and
 * locnem_samples of Accumulate_local_nematic_average (J:1009-1025). */
int j1j2c_get_locnem(void *ctx, int32_t conf, double *locspin, double *locnem, int64_t *samples);

/* Energy histogram of every slot of a conf: counts (NREPLICA x bins; bin k holds the samples of
 * J:1520-1522's histindex k+1, not yet divided by NMESS), lower edge and bin size per slot
 * (hist_en_min_t, hist_bin_size_t; any output may be NULL). */
int j1j2c_get_histogram(void *ctx, int32_t conf, double *counts, double *emin, double *binsize);

/* Recorded trace of one conf: obs (cycles x NREPLICA x 5, by slot: mag, en, strx, stry, nbar),
 * temp_of_rep (cycles x NREPLICA, by replica); *ncycles = rows written (<= trace_cycles).  The
 * per-cycle data behind cfbt / cftr (J:1397-1475) and the LOCAL lists of Process_data. */
int j1j2c_get_trace(void *ctx, int32_t conf, double *obs, int32_t *temp_of_rep, int64_t *ncycles);

/* Accepted flips per site of every slot of a conf (NREPLICA x N int32, slot-major, site order;
 * vacancies read -1 as Mark_vacancy_flipcounts sets them), counted since j1j2c_init_spins
 * (confnumflips, J:109, J:2575). */
int j1j2c_get_flip_counts(void *ctx, int32_t conf, int32_t *counts);

/* ---------------------------------------------------------------------------------------------
 * Checkpoint / resume (no reference counterpart: the reference restarts runs from scratch)
 * ------------------------------------------------------------------------------------------- */

/* Bytes of the state blob of this context. */
int j1j2c_state_size(void *ctx, int64_t *bytes);

/* Copy the whole device state into buf (at least j1j2c_state_size bytes): spins, disorder,
 * ladders, slot maps, swap counters, running sums, visit flags, last observables, cluster
 * sizes, the PT cycle counter and swap phase, and the enabled diagnostics.  Continuing a run
 * from the blob (j1j2c_load_state into a context created with the same parameters) reproduces
 * the uninterrupted run bit for bit. */
int j1j2c_save_state(void *ctx, void *buf, int64_t size);

/* Restore a blob written by j1j2c_save_state.  The context must have been created with the
 * same lattice-shape groups, couplings, precision, ptswapever, seed and conf_base
 * (J1J2C_EINVAL otherwise); the blob's diagnostics settings replace the context's. */
int j1j2c_load_state(void *ctx, const void *buf, int64_t size);

/* ---------------------------------------------------------------------------------------------
 * Results in the reference's file formats (host side; replaces the per-configuration
 * finalisation J:1542-1684, Collect_data J:2917-3207 and Write_files J:3210-3575)
 * ------------------------------------------------------------------------------------------- */

/* An accumulator of disorder averages for a run of NREPLICA temperatures temps[] (T of each slot). */
int j1j2c_results_create(void **res, const j1j2c_run_info *info, const double *temps);

/* Add one disorder configuration: its slot sums (NREPLICA records, j1j2c_get_slot_sums), occupied
 * sites (L3 - nimp), swap attempts / accepts (NREPLICA - 1 each, may be NULL), replicas that
 * visited both ladder ends, and optionally the histogram (NREPLICA x bins counts with per-slot
 * lower edge and bin size, j1j2c_get_histogram), the flip counts (NREPLICA x N,
 * j1j2c_get_flip_counts) and the random field (N). */
int j1j2c_results_add_conf(void *res, const j1j2c_slot_sums *sums, int32_t nocc,
                           const int64_t *swap_attempts, const int64_t *swap_accepts,
                           int32_t visited_both, const double *hist_counts,
                           const double *hist_min, const double *hist_bin,
                           const int32_t *flip_counts, const double *p);

/* Write cfen / cfma / cfnm / cfst / cfnd (always), cfhs (bins > 0), cfxy (write_strip),
 * cfnu (write_numflips), cfpt (PT sampler), cfph (write_phitable) into directory dir, named as
 * the reference names them (e.g. cfen00320032.dat for L = H = 32). */
int j1j2c_results_write(void *res, const char *dir);

void j1j2c_results_destroy(void *res);

/* Sweep-kernel timing accumulated under J1J2C_FLAG_PROFILE: milliseconds, launches, and the
 * attempts those launches made (occupied sites x sweeps).  Every PT cycle brackets its sweep
 * launches with its own pair of CUDA events; j1j2c_run reads them after its final
 * synchronisation, so profiling adds no host wait between the cycles of a run. */
int j1j2c_get_profile(void *ctx, double *sweep_ms, int64_t *sweep_launches, int64_t *attempts);

/* Kernel configuration the context chose: threads per CTA, sites per thread per colour phase
 * (4 = quad path, 1 = per-site path), dynamic shared memory bytes per CTA (of the first group's
 * kernel, or of the persistent launch over every group when the context uses it). */
int j1j2c_get_config(void *ctx, int32_t *block_threads, int32_t *sites_per_thread,
                     int32_t *smem_bytes);

/* ---------------------------------------------------------------------------------------------
 * Host-side model helpers (no GPU needed)
 * ------------------------------------------------------------------------------------------- */

/* make_corr_rand_3d (CR:191-386): exponential correlation of length xi on the power-of-two
 * padded periodic cube, KISS polar Gaussian noise after gkissinit(seed), Fourier filter, crop,
 * and (do_uniform) the erfcc map to [-max_value, max_value].  out[(k*n2 + j)*n1 + i] = x(i,j,k).
 * FP64 throughout. */
int j1j2c_corr_rand_3d(int32_t n1, int32_t n2, int32_t n3, double xi, int32_t seed,
                       int32_t do_uniform, double max_value, double *out);

/* Same as j1j2c_corr_rand_3d with the three 3-D transforms, the filter and the crop on the current
 * GPU (cuFFT); the white noise is drawn on the host in the reference's order and the uniform map
 * is applied on the host.  Agrees with the host form to the rounding of the transforms. */
int j1j2c_corr_rand_3d_gpu(int32_t n1, int32_t n2, int32_t n3, double xi, int32_t seed,
                           int32_t do_uniform, double max_value, double *out);

/* Setup_vacancies (J:1111-1165) after kissinit(seed): mode 0 = RAN (Bernoulli pp per site),
 * 1 = COR (anticorrelated); then bond masks with pph / ppv.  Returns the vacancy count (>= 0). */
int j1j2c_setup_vacancies(int32_t seed, int32_t L, int32_t H, double pp, double pph, double ppv,
                          int32_t mode, int8_t *occu, int8_t *jh, int8_t *jv);

/* Initialize_spin_array (J:1179-1209) after kissinit(seed), for callers that want the
 * reference's KISS-generated HOT start (then pass the result to j1j2c_init_spins). */
int j1j2c_kiss_spins(int32_t seed, int32_t L, int32_t H, int32_t start, int32_t axis, int8_t *s);

/* Temperatures of Setup_temperature_ladder (J:928-962, PT branch): split = 0 LINEAR,
 * 1 SPLIT around tmid with fraction tfrac of the intervals below it. */
int j1j2c_ladder(int32_t n, double tmin, double tmax, int32_t split, double tmid, double tfrac,
                 double *temps);

/* Exact thermal averages of a lattice with L*L*H <= 32 sites (e.g. 4 x 4 x 2) by enumerating all
 * 2^N states on the current GPU, for nbeta (1..4) inverse temperatures; the Hamiltonian is that
 * of Compute_local_field (J:2498-2541), doubled slots included.  out[b*12 + q] holds, for beta[b]:
 * q = 0 ln Z, then <e>, <e^2>, <|m|>, <m^2>, <m^4>, <|sx|>, <sx^2>, <|sy|>, <sy^2>, <nbar>,
 * <nbar^2> with per-occupied-site observables as in Measurement (J:2807-2842, J:1028-1048).
 * Allocates a small device scratch buffer.  No reference counterpart (the reference samples). */
int j1j2c_enumerate_exact(int32_t L, int32_t H, double J1h, double J1v, double J2, double J3,
                          const double *p, const int8_t *occu, const int8_t *jh,
                          const int8_t *jv, int32_t nbeta, const double *beta, double *out);

/* The same exact enumeration without any allocation, for callers that cannot allocate device
 * memory when they need it (a host framework whose memory pool already holds the whole GPU, or a
 * latency-bound loop that must not pay for an allocation).  Its scratch is a fixed device array
 * of the library: at most 512 CTAs x 4 betas x 12 partial sums plus 48 totals (about 192 KiB,
 * held by every GPU that loads the library until exit), enough for any lattice of <= 32 sites.
 * Larger requests (more than 32 sites or 4 betas) return J1J2C_EINVAL.  The first call on a
 * device looks the array's device address up (cudaGetSymbolAddress) with that device current;
 * make that first call before any stream capture.  The address is kept for the life of the
 * process, so a cudaDeviceReset between calls is not supported.  Calls share the array: calls
 * that overlap on the GPU race.  Arguments and output as j1j2c_enumerate_exact.  No counterpart
 * in the reference. */
int j1j2c_enumerate_exact_noalloc(int32_t L, int32_t H, double J1h, double J1v, double J2,
                                  double J3, const double *p, const int8_t *occu,
                                  const int8_t *jh, const int8_t *jv, int32_t nbeta,
                                  const double *beta, double *out);

/* Failure injection for tests of the error paths (process-wide, one shot): kind 1 fails the next
 * device allocation of an engine context as out of memory (J1J2C_ENOMEM from the call that made
 * it), kind 2 the next PT-cycle launch of j1j2c_run (J1J2C_ECUDA); 0 clears.  The failure is
 * reported without calling CUDA, so the device and every context stay usable.  No reference
 * counterpart (the reference stops on errors: MPI_ABORT / stop, J:443-444, J:841-925). */
int j1j2c_inject_fault(int32_t kind);

/* Library version string. */
const char *j1j2c_version(void);

#ifdef __cplusplus
}
#endif
#endif /* J1J2C_H */
