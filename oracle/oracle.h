/*
 * ORACLE — test infrastructure only.
 *
 * CPU restatement of the hot path of sim/J1J2_6tv.f90 (ShadowQFT/J1J2-public): KISS05, the
 * Metropolis sweep with the random field on the nematic variable, Measurement, the spatial mean
 * local nematic, the PT SERIAL driver and its per-slot accumulation; plus a replay of the device
 * engine's colour-ordered, Philox-keyed FP64 sweep, fixed-point energy and Philox swap.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load this library,
 * and only as the checker or the timed CPU baseline.  The product (libj1j2cuda) never links it.
 *
 * Parity pin: the disorder generator is pinned against the reference's vendored Ooura C FFT
 * (oracle/_ref, golden vectors in tests/golden/).  The Fortran program itself cannot be compiled
 * in this environment (no Fortran compiler), so the sweep/PT restatement is pinned statistically
 * against the reference's own run outputs (data/raw) and by exact enumeration.
 */
#ifndef J1J2_ORACLE_H
#define J1J2_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* lattice view for the reference-order arithmetic (site = x + L*y + L*L*z, J:539) */
typedef struct {
    int32_t L, H, N, nimp;
    double J1h, J1v, J2, J3;
    const int32_t *m;     /* 10*N neighbour table, m[k*N + i], k = 0..9 for m1..m10 (J:532-586) */
    const int8_t *occu, *jh, *jv;
    const double *p;      /* random field per site */
} or_lat;

/* number of doubles in one slot-sum record (same field order as j1j2c_slot_sums) */
#define OR_NSUM 22

/* KISS05 */
void or_kiss_init(uint32_t st[4], int32_t seed);
double or_kiss_u(uint32_t st[4]);
void or_kiss_draw(int32_t seed, int32_t n, double *out);
void or_gkiss_fill(int32_t seed, int32_t n, double *out);
double or_erfcc(double x);

/* model set-up */
void or_neighbors(int32_t L, int32_t H, int32_t *m);
int32_t or_setup_vacancies(int32_t seed, int32_t L, int32_t H, double pp, double pph, double ppv,
                           int32_t mode, const int32_t *m, int8_t *occu, int8_t *jh, int8_t *jv);
void or_init_spins(int32_t seed, int32_t L, int32_t H, int32_t start, int32_t axis, int8_t *s);
void or_ladder(int32_t n, double tmin, double tmax, int32_t split, double tmid, double tfrac,
               double *temps);

/* reference arithmetic */
double or_field_ref(const or_lat *g, const int8_t *s, int32_t i, double *n_out);
void or_measurement_ref(const or_lat *g, const int8_t *s, double out[4]);
double or_nbar_ref(const or_lat *g, const int8_t *s);
void or_metro_sweep_ref(const or_lat *g, int8_t *s, double beta, int32_t *flipcounts,
                        double obs[4], uint32_t kiss[4], int32_t rnd_order, int32_t *order);
void or_pt_serial_ref(const or_lat *g, int32_t nrep, const double *beta, int32_t ptswapever,
                      int32_t neq, int32_t nmess, int32_t irinit, int32_t iconf, int32_t start,
                      int32_t axis, double *sums, int64_t *attempts, int64_t *accepts,
                      int32_t *visitboth, int8_t *spins_out, int32_t *rep_at_temp_out);
void or_local_ref(const or_lat *g, const int8_t *s0, double beta, int32_t neq, int32_t nmess,
                  uint32_t kiss[4], double *maglist, double *enlist, double *strxlist,
                  double *strylist, double *nbarlist, int8_t *s_out);
double or_bench_pt_ref(const or_lat *g, int32_t nthreads, int32_t nrep, const double *beta,
                       int32_t ptswapever, int32_t ncycles, int32_t irinit);
double or_bench_pt_multi(const or_lat *const *gs, int32_t nlad, int32_t nthreads, int32_t nrep,
                         const double *beta, int32_t ptswapever, int32_t ncycles, int32_t irinit);

/* device-engine replay */
void or_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
double or_dexp(double x);
int64_t or_replay_sweeps(const or_lat *g, int8_t *s, double beta, uint32_t seed, uint32_t conf,
                         uint32_t rep, uint32_t sweep0, int32_t nsweeps, int32_t *flipcounts);
void or_replay_measure(const or_lat *g, const int8_t *s, int64_t ints[4], int64_t *eacc,
                       double obs[5]);
void or_replay_pt(const or_lat *g, int32_t nrep, const double *beta, int32_t ptswapever,
                  int32_t ncycles, uint32_t cycle0, uint32_t seed, uint32_t conf, int32_t measure,
                  int32_t phase0, int8_t *spins, int32_t *rep_at_temp, int32_t *temp_of_rep,
                  double *sums, int64_t *nmeas, int64_t *attempts, int64_t *accepts,
                  uint8_t *visited, double *obs_out, int32_t *flips);
int64_t or_wolff_step(const or_lat *g, int8_t *s, double beta, uint32_t seed, uint32_t conf,
                      uint32_t rep, uint32_t cycle);
void or_hot_spins_philox(int32_t L, int32_t H, uint32_t seed, uint32_t conf, uint32_t rep,
                         int8_t *s);

#ifdef __cplusplus
}
#endif
#endif
